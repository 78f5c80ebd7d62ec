"""Generate the golden fixtures in this folder from the reference itself.

Runs where the qibojit sources are available: pass the folder that holds the
``qibojit`` package (the reference's ``src`` folder) as the first argument or in
``QIBOJIT_SRC``; the GPU machine only reads the committed ``.npz`` files.  numba is not installed there, so a stand-in module with
``njit`` = identity and ``prange`` = ``range`` is placed in ``sys.modules`` first:
this is the reference CI's own ``NUMBA_DISABLE_JIT=1`` mode
(``pyproject.toml:55``), in which the kernels of
``src/qibojit/custom_operators/gates.py`` and ``ops.py`` run unchanged as Python.

The base-method arithmetic (bit position m = n-q-1, ``nstates``, ``swap_targets``,
the multi-target operand) follows ``src/qibojit/backends/cpu.py:565-635``; the case
lists follow the parametrisations of ``tests/test_gates.py`` and
``tests/test_ops.py``.  Usage: ``python tests/golden/make_golden.py <qibojit src folder>``.
"""
from __future__ import annotations

import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = None  # set by main() from the command line or QIBOJIT_SRC


def _load_reference():
    stub = types.ModuleType("numba")

    def njit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    stub.njit = njit
    stub.prange = range
    sys.modules["numba"] = stub
    mods = {}
    for name in ("gates", "ops"):
        path = os.path.join(SRC, "qibojit", "custom_operators", f"{name}.py")
        spec = importlib.util.spec_from_file_location(f"_qibojit_ref_{name}", path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mods[name] = mod
    return mods["gates"], mods["ops"]


def _rand_state(rng, n, dtype):
    x = rng.standard_normal(2**n) + 1j * rng.standard_normal(2**n)
    x /= np.linalg.norm(x)
    return x.astype(dtype)


def _rand_matrix(rng, d, dtype):
    return (rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))).astype(dtype)


def qubits_tensor(nqubits, targets, controls=()):
    q = [nqubits - t - 1 for t in targets] + [nqubits - c - 1 for c in controls]
    return np.array(sorted(q), dtype=np.int32)


def one_qubit(G, state, nqubits, target, kernel, gate, qubits):
    ncontrols = len(qubits) - 1
    m = nqubits - target - 1
    nstates = 1 << (nqubits - ncontrols - 1)
    if ncontrols:
        return getattr(G, f"multicontrol_{kernel}_kernel")(state, gate, qubits, nstates, m)
    return getattr(G, f"{kernel}_kernel")(state, gate, nstates, m)


def two_qubit(G, state, nqubits, t1, t2, kernel, gate, qubits):
    ncontrols = len(qubits) - 2
    if t1 > t2:
        swap, m1, m2 = True, nqubits - t1 - 1, nqubits - t2 - 1
    else:
        swap, m1, m2 = False, nqubits - t2 - 1, nqubits - t1 - 1
    nstates = 1 << (nqubits - 2 - ncontrols)
    if ncontrols:
        return getattr(G, f"multicontrol_{kernel}_kernel")(state, gate, qubits, nstates, m1, m2, swap)
    return getattr(G, f"{kernel}_kernel")(state, gate, nstates, m1, m2, swap)


def multi_qubit(G, state, nqubits, targets, gate, qubits):
    nstates = 1 << (nqubits - len(qubits))
    t = np.array([1 << (nqubits - q - 1) for q in targets[::-1]], dtype=np.int64)
    k = len(targets)
    kern = {3: G.apply_three_qubit_gate_kernel, 4: G.apply_four_qubit_gate_kernel,
            5: G.apply_five_qubit_gate_kernel}.get(k, G.apply_multi_qubit_gate_kernel)
    return kern(state, gate, qubits, nstates, t)


# Placement tables of tests/test_gates.py
ONE_Q = [(5, 4, []), (4, 2, []), (3, 0, []), (8, 5, []), (3, 0, [1, 2]), (4, 3, [0, 1, 2]),
         (5, 3, [1]), (5, 2, [1, 4]), (6, 3, [0, 2, 5]), (6, 3, [0, 2, 4, 5]),
         (4, 1, []), (6, 5, []), (9, 0, [8]), (9, 8, [0])]
PAULI = [(3, 0, []), (4, 3, []), (5, 2, []), (3, 1, []), (3, 0, [1]), (4, 3, [0, 1]), (5, 2, [1, 3, 4])]
ZPOW = [(3, 0, []), (3, 2, [1]), (3, 2, [0, 1]), (6, 1, [0, 2, 4])]
TWO_Q = [(5, [3, 4], []), (4, [2, 0], []), (2, [0, 1], []), (8, [6, 3], []), (3, [0, 1], [2]),
         (4, [1, 3], [0]), (5, [2, 3], [1, 4]), (5, [3, 1], [0, 2]), (6, [2, 5], [0, 1, 3, 4])]
SWAP = [(2, [0, 1], []), (3, [0, 2], []), (4, [1, 3], []), (3, [1, 2], [0]), (4, [0, 2], [1]),
        (4, [2, 3], [0]), (5, [3, 4], [1, 2]), (6, [1, 4], [0, 2, 5])]
FSIM = [(3, [0, 1], []), (4, [2, 0], []), (3, [1, 2], [0]), (4, [0, 1], [2]), (5, [0, 1], [2]),
        (5, [3, 4], [2]), (4, [0, 3], [1]), (4, [3, 2], [0]), (5, [1, 4], [2]), (6, [1, 3], [0, 4]),
        (6, [5, 0], [1, 2, 3])]
MULTI = [(3, [0, 1, 2], []), (4, [2, 1, 3], []), (5, [0, 2, 3], []), (8, [2, 6, 3], []),
         (5, [0, 2, 3, 4], []), (8, [0, 4, 2, 5, 7], []), (7, [0, 2, 4, 3, 6, 5], []),
         (8, [0, 4, 2, 3, 5, 7, 1], []), (4, [2, 1, 3], [0]), (5, [0, 2, 3], [1]),
         (8, [2, 6, 3], [4, 7]), (5, [0, 2, 3, 4], [1]), (8, [0, 4, 2, 5, 7], [1, 3]),
         (10, [0, 4, 2, 5, 9], [1, 3, 7, 8])]
COLLAPSE = [(2, [0], [1]), (2, [1], [0]), (3, [1], [1]), (4, [1, 3], [1, 0]), (5, [1, 2, 4], [0, 1, 1]),
            (10, [4, 7], [0, 0]), (11, [8, 2, 10], [1, 0, 1]), (12, [0, 1, 2, 3], [1, 0, 1, 1])]


def main():
    G, O = _load_reference()
    rng = np.random.default_rng(20261203)
    records = {}

    def put(key, **arrays):
        for name, value in arrays.items():
            records[f"{key}/{name}"] = np.asarray(value)

    idx = 0
    for dtype in ("complex128", "complex64"):
        for (n, t, c) in ONE_Q:
            for kernel in ("apply_gate", "apply_x", "apply_y", "apply_z", "apply_z_pow"):
                if kernel in ("apply_x", "apply_y", "apply_z") and (n, t, c) not in PAULI and n > 6:
                    continue
                s0 = _rand_state(rng, n, dtype)
                if kernel == "apply_gate":
                    gate = _rand_matrix(rng, 2, dtype)
                elif kernel == "apply_z_pow":
                    gate = np.asarray(np.exp(1j * rng.uniform(0, 2 * np.pi)), dtype=dtype)
                else:
                    gate = np.zeros((2, 2), dtype=dtype)
                q = qubits_tensor(n, [t], c)
                out = one_qubit(G, s0.copy(), n, t, kernel, gate, q)
                put(f"one/{idx:04d}", kernel=kernel, nqubits=n, targets=[t], controls=c, state=s0,
                    gate=gate, qubits=q, out=out)
                idx += 1
        for (n, ts, c) in TWO_Q + SWAP + FSIM:
            for kernel in ("apply_two_qubit_gate", "apply_swap", "apply_fsim"):
                s0 = _rand_state(rng, n, dtype)
                if kernel == "apply_two_qubit_gate":
                    gate = _rand_matrix(rng, 4, dtype)
                elif kernel == "apply_fsim":
                    u = _rand_matrix(rng, 2, dtype)
                    phase = np.exp(-1j * rng.uniform(0, 2 * np.pi))
                    gate = np.array([u[0, 0], u[0, 1], u[1, 0], u[1, 1], phase], dtype=dtype)
                else:
                    gate = np.zeros((4, 4), dtype=dtype)
                q = qubits_tensor(n, ts, c)
                out = two_qubit(G, s0.copy(), n, ts[0], ts[1], kernel, gate, q)
                put(f"two/{idx:04d}", kernel=kernel, nqubits=n, targets=ts, controls=c, state=s0,
                    gate=gate, qubits=q, out=out)
                idx += 1
        for (n, ts, c) in MULTI:
            s0 = _rand_state(rng, n, dtype)
            gate = _rand_matrix(rng, 2 ** len(ts), dtype)
            q = qubits_tensor(n, ts, c)
            out = multi_qubit(G, s0.copy(), n, ts, gate, q)
            put(f"multi/{idx:04d}", kernel="apply_multi_qubit_gate", nqubits=n, targets=ts, controls=c,
                state=s0, gate=gate, qubits=q, out=out)
            idx += 1
        for (n, ts, rs) in COLLAPSE:
            for normalize in (True, False):
                s0 = _rand_state(rng, n, dtype)
                q = np.array([n - t - 1 for t in reversed(sorted(ts))], dtype=np.int32)
                result = int(np.array(rs).dot(2 ** np.arange(len(rs) - 1, -1, -1)))
                fn = O.collapse_state_normalized if normalize else O.collapse_state
                out = fn(s0.copy(), q, result, n)
                put(f"collapse/{idx:04d}", nqubits=n, targets=sorted(ts), result=result,
                    normalize=normalize, state=s0, qubits=q, out=out)
                idx += 1
        s = O.initial_state_vector(np.full(16, 7, dtype=dtype))
        put(f"init/{idx:04d}", nqubits=4, out=s)
        idx += 1

    # Metropolis frequencies, ops.py:82-108 (includes the known-answer case of
    # tests/test_ops.py:236-256: uniform 16 bins, seed 1234, 4 chains, 1000 shots).
    freq_cases = [(4, 1000, 1234, 4, "uniform", "float64"), (4, 1000, 1234, 4, "uniform", "float32"),
                  (4, 1000, 1234, 1, "uniform", "float64"), (6, 5000, 42, 3, "random", "float64"),
                  (8, 20000, 7, 8, "random", "float64"), (5, 3001, 99, 5, "random", "float32"),
                  (3, 2000, 5, 2, "sparse", "float64"), (10, 10000, 123, 4, "state", "float64")]
    for (nq, nshots, seed, nthreads, kind, rt) in freq_cases:
        if kind == "uniform":
            probs = np.ones(2**nq) / 2**nq
        elif kind == "sparse":
            probs = np.zeros(2**nq)
            probs[[1, 4, 6]] = 1.0
            probs /= probs.sum()
        elif kind == "state":
            probs = np.abs(_rand_state(rng, nq, "complex128")) ** 2
        else:
            probs = rng.random(2**nq)
            probs /= probs.sum()
        probs = probs.astype(rt)
        freqs = O.measure_frequencies(np.zeros(2**nq, dtype=np.int64), probs, nshots, nq, seed, nthreads)
        put(f"freq/{idx:04d}", nqubits=nq, nshots=nshots, seed=seed, nthreads=nthreads, probs=probs,
            out=freqs)
        idx += 1

    path = os.path.join(HERE, "reference_kernels.npz")
    np.savez_compressed(path, **records)
    print(f"wrote {len(records)} arrays to {path}")


if __name__ == "__main__":
    SRC = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("QIBOJIT_SRC")
    if not SRC or not os.path.isdir(os.path.join(SRC, "qibojit")):
        sys.exit("usage: make_golden.py <folder holding the qibojit package> (or set QIBOJIT_SRC)")
    main()
