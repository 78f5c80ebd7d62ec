"""ctypes front end of the CPU oracle (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` use
this module, as the checker.  The functions keep the names and argument order of
the reference Numba kernels (``src/qibojit/custom_operators/gates.py`` and
``ops.py``) so that parity tests read like the reference's own tests; each one
mutates ``state`` in place and returns it, as the reference kernels do.

``OracleBackend`` restates the dispatch of ``NumbaBackend`` (``src/qibojit/
backends/cpu.py:433-450, 541-635``): qubit q is bit n-q-1, the ``qubits``
operand is the sorted bit positions of controls and targets, two-target gates
swap their row order when target1 > target2, and multi-target gates receive
``[1 << (n-t-1) for t in targets[::-1]]``.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

from . import build as _build

_DT = {np.dtype("complex128"): 0, np.dtype("complex64"): 1,
       np.dtype("float64"): 2, np.dtype("float32"): 3}
K_GATE, K_X, K_Y, K_Z, K_ZPOW = range(5)
K2_GATE, K2_SWAP, K2_FSIM = range(3)

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        vp, i32p, i64p = ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p
        L.oracle_one_qubit.argtypes = [ctypes.c_int, ctypes.c_int, vp, vp, i32p, ctypes.c_int,
                                       ctypes.c_int64, ctypes.c_int]
        L.oracle_two_qubit.argtypes = [ctypes.c_int, ctypes.c_int, vp, vp, i32p, ctypes.c_int,
                                       ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_multi_qubit.argtypes = [ctypes.c_int, vp, vp, i32p, ctypes.c_int, ctypes.c_int64,
                                         i64p, ctypes.c_int]
        L.oracle_initial_state.argtypes = [ctypes.c_int, vp, ctypes.c_int64]
        L.oracle_collapse_state.argtypes = [ctypes.c_int, vp, i32p, ctypes.c_int, ctypes.c_int64,
                                            ctypes.c_int, ctypes.c_int]
        L.oracle_probabilities.argtypes = [ctypes.c_int, vp, ctypes.c_int, i32p, ctypes.c_int, vp]
        L.oracle_measure_frequencies.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int64,
                                                 ctypes.c_int64, ctypes.c_uint32, ctypes.c_int, vp]
        L.oracle_mt_stream.argtypes = [ctypes.c_uint32, ctypes.c_int, ctypes.c_uint64,
                                       ctypes.c_int64, vp]
        L.oracle_multicontrol_index.argtypes = [ctypes.c_int64, i32p, ctypes.c_int]
        L.oracle_multicontrol_index.restype = ctypes.c_int64
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def max_threads() -> int:
    return lib().oracle_max_threads()


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


def _check_state(state: np.ndarray) -> int:
    if not (isinstance(state, np.ndarray) and state.flags.c_contiguous):
        raise TypeError("oracle kernels need a C-contiguous numpy array")
    return _DT[state.dtype]


def _operand(gate, dtype) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(gate, dtype=dtype).ravel())


def _qubits(qubits) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(qubits, dtype=np.int32))


def _one(kind, state, gate, qubits, nstates, m):
    dt = _check_state(state)
    g = _operand(gate if gate is not None else [0], state.dtype)
    q = _qubits(qubits if qubits is not None else [])
    rc = lib().oracle_one_qubit(dt, kind, _ptr(state), _ptr(g), _ptr(q), len(q), int(nstates), int(m))
    if rc:
        raise ValueError("oracle: unsupported dtype for this kernel")
    return state


def _two(kind, state, gate, qubits, nstates, m1, m2, swap_targets):
    dt = _check_state(state)
    g = _operand(gate if gate is not None else [0], state.dtype)
    q = _qubits(qubits if qubits is not None else [])
    rc = lib().oracle_two_qubit(dt, kind, _ptr(state), _ptr(g), _ptr(q), len(q), int(nstates),
                                int(m1), int(m2), int(bool(swap_targets)))
    if rc:
        raise ValueError("oracle: unsupported dtype")
    return state


# --- gates.py kernels (same names and argument order) -----------------------------
def apply_gate_kernel(state, gate, nstates, m):
    return _one(K_GATE, state, gate, None, nstates, m)


def multicontrol_apply_gate_kernel(state, gate, qubits, nstates, m):
    return _one(K_GATE, state, gate, qubits, nstates, m)


def apply_x_kernel(state, gate, nstates, m):
    return _one(K_X, state, None, None, nstates, m)


def multicontrol_apply_x_kernel(state, gate, qubits, nstates, m):
    return _one(K_X, state, None, qubits, nstates, m)


def apply_y_kernel(state, gate, nstates, m):
    return _one(K_Y, state, None, None, nstates, m)


def multicontrol_apply_y_kernel(state, gate, qubits, nstates, m):
    return _one(K_Y, state, None, qubits, nstates, m)


def apply_z_kernel(state, gate, nstates, m):
    return _one(K_Z, state, None, None, nstates, m)


def multicontrol_apply_z_kernel(state, gate, qubits, nstates, m):
    return _one(K_Z, state, None, qubits, nstates, m)


def apply_z_pow_kernel(state, gate, nstates, m):
    return _one(K_ZPOW, state, gate, None, nstates, m)


def multicontrol_apply_z_pow_kernel(state, gate, qubits, nstates, m):
    return _one(K_ZPOW, state, gate, qubits, nstates, m)


def apply_two_qubit_gate_kernel(state, gate, nstates, m1, m2, swap_targets=False):
    return _two(K2_GATE, state, gate, None, nstates, m1, m2, swap_targets)


def multicontrol_apply_two_qubit_gate_kernel(state, gate, qubits, nstates, m1, m2, swap_targets=False):
    return _two(K2_GATE, state, gate, qubits, nstates, m1, m2, swap_targets)


def apply_swap_kernel(state, gate, nstates, m1, m2, swap_targets=False):
    return _two(K2_SWAP, state, None, None, nstates, m1, m2, swap_targets)


def multicontrol_apply_swap_kernel(state, gate, qubits, nstates, m1, m2, swap_targets=False):
    return _two(K2_SWAP, state, None, qubits, nstates, m1, m2, swap_targets)


def apply_fsim_kernel(state, gate, nstates, m1, m2, swap_targets=False):
    return _two(K2_FSIM, state, gate, None, nstates, m1, m2, swap_targets)


def multicontrol_apply_fsim_kernel(state, gate, qubits, nstates, m1, m2, swap_targets=False):
    return _two(K2_FSIM, state, gate, qubits, nstates, m1, m2, swap_targets)


def apply_multi_qubit_gate_kernel(state, gate, qubits, nstates, targets):
    dt = _check_state(state)
    g = _operand(gate, state.dtype)
    q = _qubits(qubits)
    t = np.ascontiguousarray(np.asarray(targets, dtype=np.int64))
    if g.size != (1 << (2 * len(t))):
        raise ValueError("gate size does not match the number of targets")
    lib().oracle_multi_qubit(dt, _ptr(state), _ptr(g), _ptr(q), len(q), int(nstates), _ptr(t), len(t))
    return state


apply_three_qubit_gate_kernel = apply_multi_qubit_gate_kernel
apply_four_qubit_gate_kernel = apply_multi_qubit_gate_kernel
apply_five_qubit_gate_kernel = apply_multi_qubit_gate_kernel


def multicontrol_index(g, qubits):
    q = _qubits(qubits)
    return lib().oracle_multicontrol_index(int(g), _ptr(q), len(q))


# --- ops.py -------------------------------------------------------------------------
def initial_state_vector(state):
    dt = _check_state(state)
    lib().oracle_initial_state(dt, _ptr(state), state.size)
    return state


def collapse_state(state, qubits, result, nqubits):
    dt = _check_state(state)
    q = _qubits(qubits)
    lib().oracle_collapse_state(dt, _ptr(state), _ptr(q), len(q), int(result), int(nqubits), 0)
    return state


def collapse_state_normalized(state, qubits, result, nqubits):
    dt = _check_state(state)
    q = _qubits(qubits)
    lib().oracle_collapse_state(dt, _ptr(state), _ptr(q), len(q), int(result), int(nqubits), 1)
    return state


def measure_frequencies(frequencies, probs, nshots, nqubits, seed, nthreads):
    """ops.py:82-108.  Accumulates into ``frequencies`` (any integer dtype) and returns it."""
    p = np.ascontiguousarray(probs)
    if p.dtype == np.float64:
        rt = 0
    elif p.dtype == np.float32:
        rt = 1
    else:
        raise TypeError("probs must be float32 or float64")
    f64 = np.zeros(frequencies.shape[0], dtype=np.int64)
    rc = lib().oracle_measure_frequencies(_ptr(f64), _ptr(p), rt, frequencies.shape[0], int(nshots),
                                          int(seed) & 0xFFFFFFFF, int(nthreads), None)
    if rc:
        raise ValueError("oracle measure_frequencies: bad arguments or out of memory")
    frequencies += f64.astype(frequencies.dtype)
    return frequencies


def chain_seeds(seed: int, nthreads: int) -> np.ndarray:
    """The per-chain seeds ops.py:92-93 draws (np.random.seed(seed); randint(0, 1e8) each)."""
    out = np.zeros(nthreads, dtype=np.uint32)
    f = np.zeros(1, dtype=np.int64)
    p = np.ones(1, dtype=np.float64)
    lib().oracle_measure_frequencies(_ptr(f), _ptr(p), 0, 1, 0, int(seed) & 0xFFFFFFFF, int(nthreads),
                                     _ptr(out))
    return out


def mt_stream(seed: int, kind: str, count: int, high: int = 0) -> np.ndarray:
    code = {"word": 0, "randint": 1, "random": 2}[kind]
    out = np.zeros(count, dtype=np.float64)
    lib().oracle_mt_stream(int(seed) & 0xFFFFFFFF, code, int(high), int(count), _ptr(out))
    return out


def sample_shots(probs: np.ndarray, uniforms: np.ndarray) -> np.ndarray:
    """Direct sampling as the reference's branch below SHOT_METROPOLIS_THRESHOLD
    (``cpu.py:384-385``) reaches it: qibo's ``Backend.sample_shots`` is
    ``numpy.random.choice(N, nshots, p=probs)``, whose legacy algorithm normalises
    ``cdf = cumsum(p) / cdf[-1]`` in FP64, draws one ``random_sample`` per shot and
    returns ``cdf.searchsorted(u, side="right")``.  The caller passes those uniforms."""
    cdf = np.cumsum(np.asarray(probs, dtype=np.float64))
    cdf /= cdf[-1]
    return np.searchsorted(cdf, np.asarray(uniforms, dtype=np.float64), side="right").astype(np.int64)


def probabilities(state: np.ndarray, qubits: Sequence[int], nqubits: int) -> np.ndarray:
    """|psi|^2 marginalised on ``qubits`` (qubit indices, qubits[0] most significant)."""
    dt = _check_state(state)
    q = _qubits(list(qubits))
    out = np.zeros(1 << len(q), dtype=np.float64)
    lib().oracle_probabilities(dt, _ptr(state), int(nqubits), _ptr(q), len(q), _ptr(out))
    return out


# --- NumbaBackend dispatch (cpu.py:433-450, 541-635) ---------------------------------
class OracleBackend:
    """The reference's ``_one/_two/_multi_qubit_base`` and collapse dispatch on numpy arrays."""

    platform = "oracle"

    def __init__(self, nthreads: Optional[int] = None):
        if nthreads:
            set_threads(nthreads)

    @staticmethod
    def qubits_tensor(nqubits, targets, controls=()):
        q = [nqubits - t - 1 for t in targets] + [nqubits - c - 1 for c in controls]
        return np.array(sorted(q), dtype=np.int32)

    def _one_qubit_base(self, state, nqubits, target, kernel, gate, qubits):
        ncontrols = len(qubits) - 1 if qubits is not None else 0
        m = nqubits - target - 1
        nstates = 1 << (nqubits - ncontrols - 1)
        if ncontrols:
            return globals()[f"multicontrol_{kernel}_kernel"](state, gate, qubits, nstates, m)
        return globals()[f"{kernel}_kernel"](state, gate, nstates, m)

    def _two_qubit_base(self, state, nqubits, target1, target2, kernel, gate, qubits):
        ncontrols = len(qubits) - 2 if qubits is not None else 0
        if target1 > target2:
            swap_targets = True
            m1, m2 = nqubits - target1 - 1, nqubits - target2 - 1
        else:
            swap_targets = False
            m1, m2 = nqubits - target2 - 1, nqubits - target1 - 1
        nstates = 1 << (nqubits - 2 - ncontrols)
        if ncontrols:
            return globals()[f"multicontrol_{kernel}_kernel"](state, gate, qubits, nstates, m1, m2,
                                                               swap_targets)
        return globals()[f"{kernel}_kernel"](state, gate, nstates, m1, m2, swap_targets)

    def _multi_qubit_base(self, state, nqubits, targets, gate, qubits):
        if qubits is None:
            qubits = np.array(sorted(nqubits - q - 1 for q in targets), dtype=np.int32)
        nstates = 1 << (nqubits - len(qubits))
        t = np.array([1 << (nqubits - t - 1) for t in targets[::-1]], dtype=np.int64)
        return apply_multi_qubit_gate_kernel(state, gate, qubits, nstates, t)

    def collapse_state(self, state, qubits, shot, nqubits, normalize=True):
        q = np.array([nqubits - q - 1 for q in reversed(qubits)], dtype=np.int32)
        shot = int(np.asarray(shot).ravel()[0])
        if normalize:
            return collapse_state_normalized(state, q, shot, nqubits)
        return collapse_state(state, q, shot, nqubits)

    def zero_state(self, nqubits, dtype="complex128"):
        return initial_state_vector(np.empty(1 << nqubits, dtype=dtype))


# --- density matrices ---------------------------------------------------------------
def apply_gate_density_matrix(backend: OracleBackend, rho: np.ndarray, nqubits: int, targets, controls,
                              kernel: str, gate) -> np.ndarray:
    """rho -> U rho U^dagger on the 2n-qubit vector of the row-major rho, as
    ``_apply_gate_density_matrix`` / ``_apply_ygate_density_matrix`` (cpu.py:452-517):
    the gate's kernel with ``qubits + n`` on the row qubits, then with conj(gate) and
    ``qubits`` on the column qubits ``t + n``.  Y and CY run ``apply_y`` on the rows and
    ``apply_gate`` with conj(Y) on the columns.  ``kernel`` is the one- or two-target
    kernel name, or "multi" for ``_multi_qubit_base``."""
    flat = rho.reshape(-1)
    qubits = backend.qubits_tensor(nqubits, targets, controls)
    qubits_dm = qubits + nqubits
    targets_dm = [t + nqubits for t in targets]
    n2 = 2 * nqubits
    conj = np.conj(gate) if isinstance(gate, np.ndarray) or np.iscomplexobj(gate) else gate
    if kernel == "apply_y":
        backend._one_qubit_base(flat, n2, targets[0], "apply_y", gate, qubits_dm)
        backend._one_qubit_base(flat, n2, targets_dm[0], "apply_gate", np.conj(gate), qubits)
    elif kernel == "multi":
        backend._multi_qubit_base(flat, n2, list(targets), gate, qubits_dm)
        backend._multi_qubit_base(flat, n2, targets_dm, conj, qubits)
    elif len(targets) == 1:
        backend._one_qubit_base(flat, n2, targets[0], kernel, gate, qubits_dm)
        backend._one_qubit_base(flat, n2, targets_dm[0], kernel, conj, qubits)
    else:
        backend._two_qubit_base(flat, n2, targets[0], targets[1], kernel, gate, qubits_dm)
        backend._two_qubit_base(flat, n2, targets_dm[0], targets_dm[1], kernel, conj, qubits)
    return rho


def apply_channel_density_matrix(rho: np.ndarray, coefficients: Sequence[float], branches) -> np.ndarray:
    """``_apply_channel_density_matrix`` (cpu.py:400-415): (1 - sum c) rho + sum_k c_k
    U_k rho U_k^dagger.  ``branches[k]`` applies U_k to a density matrix in place; every
    branch starts from a copy of rho (the reference undoes unitary branches with the
    inverse gate instead, which agrees to rounding)."""
    new = (1 - float(sum(coefficients))) * rho
    for c, apply in zip(coefficients, branches):
        work = rho.copy()
        apply(work)
        new += float(c) * work
    return new


def density_probabilities(rho: np.ndarray, qubits: Sequence[int], nqubits: int) -> np.ndarray:
    """Re diag(rho) marginalised on ``qubits``, ordered as given (qubits[0] the most
    significant output bit), summed in FP64: the density-matrix branch of qibo's
    ``calculate_probabilities`` (a third-party method, restated from its definition)."""
    d = np.real(np.diagonal(np.asarray(rho).reshape(1 << nqubits, 1 << nqubits))).astype(np.float64)
    d = d.reshape((2,) * nqubits)
    rest = tuple(q for q in range(nqubits) if q not in qubits)
    marg = d.sum(axis=rest) if rest else d
    kept = [q for q in range(nqubits) if q in qubits]  # axes left, ascending
    marg = np.transpose(marg, [kept.index(q) for q in qubits])
    return np.ascontiguousarray(marg).reshape(-1)


def collapse_density_matrix(rho: np.ndarray, qubits: Sequence[int], shot: int, nqubits: int,
                            normalize: bool = True) -> np.ndarray:
    """P rho P (/ tr(P rho P)) in place, P projecting ``qubits`` onto the bits of ``shot``
    (qubits[0] its most significant bit): qibo's density-matrix collapse, restated."""
    dim = 1 << nqubits
    m = np.asarray(rho).reshape(dim, dim)
    idx = np.arange(dim)
    keep = np.ones(dim, dtype=bool)
    k = len(qubits)
    for j, q in enumerate(qubits):
        bit = (shot >> (k - 1 - j)) & 1
        keep &= ((idx >> (nqubits - 1 - q)) & 1) == bit
    p = float(np.sum(np.real(np.diagonal(m))[keep], dtype=np.float64))
    m[~keep, :] = 0
    m[:, ~keep] = 0
    if normalize:
        with np.errstate(divide="ignore", invalid="ignore"):
            m *= np.float64(1.0) / np.float64(p)
    return rho
